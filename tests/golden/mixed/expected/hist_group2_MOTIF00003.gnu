set output "hist_group2_MOTIF00003.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-20.6011:7.85821]
set yrange [0:235018]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group2_MOTIF00003.dat" using 1:2 title 'MOTIF00003 (group2)' with boxes
