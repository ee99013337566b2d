set output "hist_group1_MOTIF00008.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-32.1444:8.94594]
set yrange [0:122337]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group1_MOTIF00008.dat" using 1:2 title 'MOTIF00008 (group1)' with boxes
