set output "hist_group2_MOTIF00009.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-36.9569:11.2183]
set yrange [0:121003]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group2_MOTIF00009.dat" using 1:2 title 'MOTIF00009 (group2)' with boxes
