set output "hist_group1_MOTIF00009.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-37.0943:9.54242]
set yrange [0:108632]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group1_MOTIF00009.dat" using 1:2 title 'MOTIF00009 (group1)' with boxes
